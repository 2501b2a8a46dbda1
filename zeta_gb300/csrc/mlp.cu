/*
 * mlp.cu -- the learned move-ordering network on Blackwell tensor cores.
 *
 * Network (the project's addition; the reference orders moves by hand,
 * zeta.cl:2039-2110): 768 one-hot inputs (12 piece kinds x 64 squares,
 * from the side to move, board mirrored for black) -> 512 ReLU -> 256 ReLU
 * -> 128 = (q_from, q_to), and a move's score is
 * q_from . E_from[from] + q_to . E_to[to] with learned 64-wide square
 * embeddings.  Training minimises the softmax cross-entropy of the legal
 * moves against the best move of a plain search.
 *
 * Every matrix product -- forward, input gradients, weight gradients -- is
 * one kernel, k_gemm: C[M x N] = A[M x K] . B[N x K]^T with both operands
 * K-major BF16 (or FP8 E4M3 for inference), FP32 accumulation in tensor
 * memory.  A CTA owns a 128-row by BN-column output tile: its threads
 * stage 64-element (BF16) or 128-element (FP8) K slices of A and B into
 * 128-byte-swizzled shared memory, one thread issues the tcgen05.mma
 * instructions and commits them to an mbarrier, and after the K loop the
 * four warps read their 32 accumulator lanes back with tcgen05.ld and
 * apply the epilogue (bias, ReLU, FP32 / BF16 / transposed BF16 stores).
 * Every wait is bounded; a timeout sets an error word and the kernel
 * still frees its tensor memory.
 */
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_bf16.h>
#include <cuda_fp8.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <vector>

#include "context.cuh"
#include "tc.cuh"

namespace zeta {

namespace {

typedef __nv_bfloat16 bf16;
constexpr uint32_t kWaitTries = 1u << 22;
constexpr uint32_t MST_TIMEOUT = 1u;

struct GemmArgs {
  const void *A;      /* M x K, K-major */
  const void *B;      /* N x K, K-major */
  int M, N, K;
  const float *bias;  /* N, or null */
  int relu;
  float *Cf;          /* M x N fp32 (ldc = N), or null */
  bf16 *Cb;           /* M x N bf16, or null */
  bf16 *Ct;           /* N x M bf16 (transposed), or null */
  float scale;        /* multiplies the accumulator (FP8 dequantisation) */
  uint32_t *err;
  const bf16 *mask;   /* M x N: zero where mask <= 0 (ReLU derivative), or null */
  const unsigned *amaxA, *amaxB; /* FP8: per-tensor max |x| (float bits); scale *= amaxA*amaxB/448^2 */
};

/* The product C[M x N] = A[M x K] . B[N x K]^T of one 128 x BN output
 * tile (a K range of it when split-K), 128 threads:
 *   thread 0   TMA producer: 128-byte-wide K slices of A and B into a ring
 *              of `stages` shared-memory slots (128-byte swizzle, the
 *              layout the MMA descriptors expect), one mbarrier per slot
 *              counting the bytes in flight;
 *   thread 32  MMA issuer: four tcgen05.mma per slot into the FP32
 *              accumulator in tensor memory, then tcgen05.commit on the
 *              slot's "empty" barrier so the producer can refill it, and
 *              a final commit on `done`;
 *   all warps  epilogue: warp w reads accumulator lanes 32w..32w+31 with
 *              tcgen05.ld and applies scale, bias, ReLU, ReLU mask and the
 *              FP32 / BF16 / transposed BF16 stores (atomic FP32 adds when
 *              the K range is split across CTAs).
 * Loads of slot s+stages overlap the MMAs of slot s.  Every wait is
 * bounded: a timeout sets an error word, the producer's copies still in
 * flight are awaited (bounded), tensor memory is freed. */
constexpr int kMaxStages = 8;

/* Epilogue of one 128 x BN accumulator: the calling warp's 32 TMEM lanes
 * (tacc addresses lane 0 of them and the accumulator's first column) are
 * rows row..row of C (one row per thread); scale, bias, ReLU, ReLU mask,
 * then the FP32 / BF16 / transposed BF16 stores (atomic FP32 adds when the
 * K range was split across CTAs). */
template <int BN>
__device__ __forceinline__ void gemm_epilogue(const GemmArgs &g, uint32_t tacc, int row, int n0, float scale,
                                              bool split) {
#pragma unroll 1
  for (int c0 = 0; c0 < BN; c0 += 16) {
    float v[16];
    tc::tmem_ld16(tacc + (uint32_t)c0, v);
    const int cb = n0 + c0;
    if (row >= g.M || cb >= g.N) continue;
    const bool whole = cb + 16 <= g.N;
#pragma unroll
    for (int j = 0; j < 16; j++) {
      float x = v[j] * scale;
      if (g.bias && cb + j < g.N) x += g.bias[cb + j];
      if (g.relu) x = fmaxf(x, 0.f);
      v[j] = x;
    }
    if (g.mask) {
      const bf16 *mk = g.mask + (size_t)row * g.N + cb;
#pragma unroll
      for (int j = 0; j < 16; j++)
        if (cb + j < g.N && !(__bfloat162float(mk[j]) > 0.f)) v[j] = 0.f;
    }
    if (g.Cf) {
      float *cp = g.Cf + (size_t)row * g.N + cb;
      if (split) {
#pragma unroll
        for (int j = 0; j < 16; j++)
          if (cb + j < g.N) atomicAdd(cp + j, v[j]);
      } else if (whole && ((uintptr_t)cp & 15) == 0) {
#pragma unroll
        for (int j = 0; j < 16; j += 4) *(float4 *)(cp + j) = make_float4(v[j], v[j + 1], v[j + 2], v[j + 3]);
      } else {
#pragma unroll
        for (int j = 0; j < 16; j++)
          if (cb + j < g.N) cp[j] = v[j];
      }
    }
    if (g.Cb) {
      bf16 *cp = g.Cb + (size_t)row * g.N + cb;
      if (whole && ((uintptr_t)cp & 15) == 0) {
        __align__(16) bf16 h[16];
#pragma unroll
        for (int j = 0; j < 16; j++) h[j] = __float2bfloat16(v[j]);
        *(uint4 *)cp = *(const uint4 *)h;
        *(uint4 *)(cp + 8) = *(const uint4 *)(h + 8);
      } else {
#pragma unroll
        for (int j = 0; j < 16; j++)
          if (cb + j < g.N) cp[j] = __float2bfloat16(v[j]);
      }
    }
    if (g.Ct) {
#pragma unroll
      for (int j = 0; j < 16; j++)
        if (cb + j < g.N) g.Ct[(size_t)(cb + j) * g.M + row] = __float2bfloat16(v[j]);
    }
  }
}

__device__ __forceinline__ float gemm_scale(const GemmArgs &g) {
  float scale = g.scale;
  if (g.amaxA && g.amaxB) scale *= (__uint_as_float(*g.amaxA) / 448.f) * (__uint_as_float(*g.amaxB) / 448.f);
  return scale;
}

template <int BN, bool FP8>
__global__ void __launch_bounds__(128, 1)
    k_gemm(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB, GemmArgs g,
           int kb_per_split, int stages) {
  extern __shared__ uint8_t smem_raw[];
  uint8_t *base = (uint8_t *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  constexpr uint32_t A_BYTES = 128 * 128, B_BYTES = BN * 128, STAGE = A_BYTES + B_BYTES;
  __shared__ uint64_t full[kMaxStages], empty[kMaxStages], done;
  __shared__ uint32_t s_taddr;
  __shared__ int s_fail, s_issued;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int m0 = blockIdx.x * 128, n0 = blockIdx.y * BN;
  constexpr int EK = FP8 ? 128 : 64; /* K elements per 128-byte row */
  constexpr uint32_t IDESC = FP8 ? tc::idesc_f8(128, BN) : tc::idesc_f16(128, BN, 1);
  const int nkb = g.K / EK;
  const int kb0 = blockIdx.z * kb_per_split;
  const int cnt = min(nkb, kb0 + kb_per_split) - kb0;

  if (warp == 0) tc::tmem_alloc(&s_taddr, BN);
  if (tid == 0) {
    for (int s = 0; s < stages; s++) {
      tc::mbar_init(&full[s], 1);
      tc::mbar_init(&empty[s], 1);
    }
    tc::mbar_init(&done, 1);
    s_fail = 0;
    s_issued = 0;
    tc::prefetch_tmap(&tmA);
    tc::prefetch_tmap(&tmB);
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t taddr = s_taddr;

  if (tid == 0) {
    /* producer */
    int i = 0;
    for (; i < cnt; i++) {
      const int s = i % stages;
      if (i >= stages && !tc::mbar_wait(&empty[s], ((i / stages) - 1) & 1, kWaitTries)) {
        s_fail = 1;
        break;
      }
      uint8_t *sa = base + (size_t)s * STAGE;
      tc::mbar_arrive_expect_tx(&full[s], STAGE);
      tc::tma_load_2d(sa, &tmA, (kb0 + i) * EK, m0, &full[s]);
      tc::tma_load_2d(sa + A_BYTES, &tmB, (kb0 + i) * EK, n0, &full[s]);
    }
    s_issued = i;
  } else if (tid == 32) {
    /* MMA issuer */
    for (int i = 0; i < cnt; i++) {
      const int s = i % stages;
      if (!tc::mbar_wait(&full[s], (i / stages) & 1, kWaitTries)) {
        s_fail = 1;
        break;
      }
      tc::fence_after_sync();
      const uint32_t a0 = tc::smem_u32(base + (size_t)s * STAGE), b0 = a0 + A_BYTES;
#pragma unroll
      for (int j = 0; j < 4; j++) {
        const uint64_t ad = tc::smem_desc_sw128(a0 + 32 * j), bd = tc::smem_desc_sw128(b0 + 32 * j);
        if (FP8) tc::mma_f8(taddr, ad, bd, IDESC, (i > 0 || j > 0) ? 1u : 0u);
        else tc::mma_f16(taddr, ad, bd, IDESC, (i > 0 || j > 0) ? 1u : 0u);
      }
      tc::mma_commit(&empty[s]);
    }
    tc::mma_commit(&done); /* arrives when every MMA above has completed */
  }
  const bool finished = tc::mbar_wait(&done, 0, kWaitTries);
  __syncthreads();
  tc::fence_after_sync();
  if (finished && !s_fail) {
    gemm_epilogue<BN>(g, taddr + ((uint32_t)(warp * 32) << 16), m0 + warp * 32 + lane, n0, gemm_scale(g),
                      gridDim.z > 1);
  } else {
    if (tid == 0) {
      atomicOr(g.err, MST_TIMEOUT);
      /* copies still in flight land before the memory goes away */
      const int issued = s_issued;
      for (int i = max(0, issued - stages); i < issued; i++)
        tc::mbar_wait(&full[i % stages], (i / stages) & 1, kWaitTries);
    }
    if (tid == 32) tc::mbar_wait(&done, 0, kWaitTries);
  }
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) tc::tmem_free(taddr, BN);
}

/* The same product as a persistent kernel: one CTA per SM walks the
 * output tiles t = blockIdx.x, blockIdx.x + gridDim.x, ... (tile t is rows
 * 128 (t / nt), columns BN (t % nt), so neighbouring CTAs share their A
 * rows in L2), 192 threads:
 *   warp 0, lane 0  TMA producer: K slices of every tile in turn into a
 *                   ring of `stages` slots that runs on across tiles;
 *   warp 1, lane 0  MMA issuer: tile j into tensor-memory accumulator
 *                   j & 1 (two accumulators of BN columns), then
 *                   tcgen05.commit on that accumulator's "full" barrier;
 *   warps 2-5       epilogue: warp w reads TMEM lanes 32 (w % 4) .. + 31
 *                   of the finished accumulator, stores the rows and
 *                   releases the accumulator ("empty" barrier, one arrival
 *                   per warp).
 * So the epilogue of tile j runs under the MMAs of tile j + 1 and the
 * loads of the tiles after it.  Every wait is bounded; a timeout sets an
 * error word, every role stops, the producer's copies still in flight and
 * the issued MMAs are awaited (bounded), and tensor memory is freed.  The
 * launch asks for enough shared memory that two CTAs never share an SM,
 * so the 2 x BN-column allocation never waits for another CTA. */
constexpr int kPersistThreads = 192;
constexpr int kPersistMaxSlices = 32; /* automatic choice: persistent up to this many K slices per tile */

template <int BN, bool FP8>
__global__ void __launch_bounds__(kPersistThreads, 1)
    k_gemm_persist(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB, GemmArgs g,
                   int stages) {
  extern __shared__ uint8_t smem_raw[];
  uint8_t *base = (uint8_t *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  constexpr uint32_t A_BYTES = 128 * 128, B_BYTES = BN * 128, STAGE = A_BYTES + B_BYTES;
  __shared__ uint64_t full[kMaxStages], empty[kMaxStages], acc_full[2], acc_empty[2], done;
  __shared__ uint32_t s_taddr;
  __shared__ int s_fail;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  constexpr int EK = FP8 ? 128 : 64; /* K elements per 128-byte row */
  constexpr uint32_t IDESC = FP8 ? tc::idesc_f8(128, BN) : tc::idesc_f16(128, BN, 1);
  const int nkb = g.K / EK;
  const int nt = (g.N + BN - 1) / BN;
  const int ntiles = ((g.M + 127) / 128) * nt;

  if (warp == 0) tc::tmem_alloc(&s_taddr, 2 * BN);
  if (tid == 32) {
    for (int i = 0; i < stages; i++) {
      tc::mbar_init(&full[i], 1);
      tc::mbar_init(&empty[i], 1);
    }
    for (int a = 0; a < 2; a++) {
      tc::mbar_init(&acc_full[a], 1);
      tc::mbar_init(&acc_empty[a], 4);
    }
    tc::mbar_init(&done, 1);
    s_fail = 0;
    tc::prefetch_tmap(&tmA);
    tc::prefetch_tmap(&tmB);
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t taddr = s_taddr;
  volatile int *fail = &s_fail;

  if (warp == 0) {
    if (lane == 0) {
      /* producer */
      uint32_t it = 0;
      bool ok = true;
      for (int t = blockIdx.x; ok && t < ntiles; t += gridDim.x) {
        const int m0 = (t / nt) * 128, n0 = (t % nt) * BN;
        for (int kb = 0; kb < nkb; kb++) {
          const uint32_t sl = it % (uint32_t)stages, use = it / (uint32_t)stages;
          if ((use > 0 && !tc::mbar_wait(&empty[sl], (use - 1) & 1, kWaitTries)) || *fail) {
            ok = false;
            break;
          }
          uint8_t *sa = base + (size_t)sl * STAGE;
          tc::mbar_arrive_expect_tx(&full[sl], STAGE);
          tc::tma_load_2d(sa, &tmA, kb * EK, m0, &full[sl]);
          tc::tma_load_2d(sa + A_BYTES, &tmB, kb * EK, n0, &full[sl]);
          it++;
        }
      }
      if (!ok) {
        *fail = 1;
        /* copies still in flight land before the memory goes away */
        for (uint32_t i = it > (uint32_t)stages ? it - (uint32_t)stages : 0u; i < it; i++)
          tc::mbar_wait(&full[i % (uint32_t)stages], (i / (uint32_t)stages) & 1, kWaitTries);
      }
    }
  } else if (warp == 1) {
    if (lane == 0) {
      /* MMA issuer */
      uint32_t it = 0;
      bool ok = true;
      int j = 0;
      for (int t = blockIdx.x; ok && t < ntiles; t += gridDim.x, j++) {
        const int a = j & 1;
        if (j >= 2 && !tc::mbar_wait(&acc_empty[a], ((j >> 1) - 1) & 1, kWaitTries)) {
          ok = false;
          break;
        }
        tc::fence_after_sync();
        const uint32_t tacc = taddr + (uint32_t)(a * BN);
        for (int kb = 0; kb < nkb; kb++) {
          const uint32_t sl = it % (uint32_t)stages;
          if (!tc::mbar_wait(&full[sl], (it / (uint32_t)stages) & 1, kWaitTries) || *fail) {
            ok = false;
            break;
          }
          tc::fence_after_sync();
          const uint32_t a0 = tc::smem_u32(base + (size_t)sl * STAGE), b0 = a0 + A_BYTES;
#pragma unroll
          for (int k = 0; k < 4; k++) {
            const uint64_t ad = tc::smem_desc_sw128(a0 + 32 * k), bd = tc::smem_desc_sw128(b0 + 32 * k);
            if (FP8) tc::mma_f8(tacc, ad, bd, IDESC, (kb > 0 || k > 0) ? 1u : 0u);
            else tc::mma_f16(tacc, ad, bd, IDESC, (kb > 0 || k > 0) ? 1u : 0u);
          }
          tc::mma_commit(&empty[sl]);
          it++;
        }
        if (!ok) break;
        tc::mma_commit(&acc_full[a]); /* arrives when the tile's MMAs have completed */
      }
      if (!ok) *fail = 1;
      tc::mma_commit(&done);
      tc::mbar_wait(&done, 0, kWaitTries); /* every MMA issued above has completed */
    }
  } else {
    /* epilogue: TMEM lanes 32 q .. 32 q + 31 are rows 32 q .. of the tile */
    const int q = warp & 3;
    const float scale = gemm_scale(g);
    int j = 0;
    for (int t = blockIdx.x; t < ntiles; t += gridDim.x, j++) {
      const int a = j & 1;
      const bool got = tc::mbar_wait(&acc_full[a], (j >> 1) & 1, kWaitTries);
      /* warp-uniform decision: tcgen05.ld needs the whole warp */
      if (!__all_sync(0xFFFFFFFFu, got) || __shfl_sync(0xFFFFFFFFu, *fail, 0)) {
        if (lane == 0) *fail = 1;
        break;
      }
      tc::fence_after_sync();
      gemm_epilogue<BN>(g, taddr + ((uint32_t)(q * 32) << 16) + (uint32_t)(a * BN), (t / nt) * 128 + q * 32 + lane,
                        (t % nt) * BN, scale, false);
      tc::fence_before_sync();
      __syncwarp();
      if (lane == 0) tc::mbar_arrive(&acc_empty[a]);
    }
  }
  tc::fence_before_sync();
  __syncthreads();
  if (tid == 0 && *fail) atomicOr(g.err, MST_TIMEOUT);
  if (warp == 0) tc::tmem_free(taddr, 2 * BN);
}

/* driver's tensor-map encoder, looked up once through the runtime */
PFN_cuTensorMapEncodeTiled_v12000 tmap_encoder() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  if (!fn) {
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = (PFN_cuTensorMapEncodeTiled_v12000)p;
  }
  return fn;
}

/* a K-major operand (rows x K) as a tensor map of 128-byte-wide boxes of
 * box_rows rows, 128-byte swizzle; rows beyond the operand read as zero */
int make_tmap(CUtensorMap *m, const void *ptr, uint64_t rows, uint64_t K, int esz, uint32_t box_rows) {
  PFN_cuTensorMapEncodeTiled_v12000 enc = tmap_encoder();
  if (!enc) return set_error(ZETA_ERR_CUDA, "cuTensorMapEncodeTiled is not available");
  if (((uintptr_t)ptr & 15) || ((K * esz) & 15)) return set_error(ZETA_ERR_ARG, "gemm operand not 16-byte aligned");
  cuuint64_t dims[2] = {(cuuint64_t)K, (cuuint64_t)rows};
  cuuint64_t strides[1] = {(cuuint64_t)K * esz};
  cuuint32_t box[2] = {(cuuint32_t)(128 / esz), box_rows};
  cuuint32_t estr[2] = {1, 1};
  CUresult r = enc(m, esz == 2 ? CU_TENSOR_MAP_DATA_TYPE_BFLOAT16 : CU_TENSOR_MAP_DATA_TYPE_UINT8, 2,
                   const_cast<void *>(ptr), dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                   CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return set_error(ZETA_ERR_CUDA, "cuTensorMapEncodeTiled failed (%d)", (int)r);
  return ZETA_OK;
}

constexpr size_t gemm_stage_bytes(int BN) { return (size_t)(128 + BN) * 128; }

/* kernel choice: 0 = automatic (the persistent kernel for short K -- up to
 * kPersistMaxSlices K slices per tile, the network's shapes, where the
 * epilogue is a large share of a tile's time -- else the per-tile kernel,
 * its ring sized for 2 CTAs per SM, or 1 for split-K launches);
 * 1 or 2 = the per-tile kernel with its ring sized for 1 or 2 resident
 * CTAs per SM; 3 = the persistent kernel (split-K launches keep the
 * per-tile one) */
int g_gemm_ctas_per_sm = 0;

}  // namespace

int gemm_set_ctas_per_sm(int c) {
  if (c < 0 || c > 3)
    return set_error(ZETA_ERR_ARG, "gemm: 0 (auto), 1 or 2 (per-tile kernel, CTAs per SM) or 3 (persistent)");
  g_gemm_ctas_per_sm = c;
  return ZETA_OK;
}

/* C = A . B^T (+bias, relu) on the tensor cores; operands K-major, K a
 * multiple of 64 (BF16) or 128 (FP8), N a multiple of 16.  When only an
 * FP32 output is written and the output is small next to K (weight
 * gradients), the K range is split over CTAs that add their partial
 * products atomically; the caller zeroes C first (accumulate = 1). */
int gemm_launch(const GemmArgs &g, bool fp8, cudaStream_t s, int accumulate = 0) {
  if (g.M <= 0 || g.N <= 0 || g.K <= 0 || (g.K % (fp8 ? 128 : 64)) || (g.N % 16))
    return set_error(ZETA_ERR_ARG, "gemm: M %d N %d K %d not supported", g.M, g.N, g.K);
  const int BN = g.N >= 256 ? 256 : (g.N > 64 ? 128 : 64);
  const int esz = fp8 ? 1 : 2;
  CUtensorMap ta, tb;
  int rc = make_tmap(&ta, g.A, (uint64_t)g.M, (uint64_t)g.K, esz, 128);
  if (rc) return rc;
  rc = make_tmap(&tb, g.B, (uint64_t)g.N, (uint64_t)g.K, esz, (uint32_t)BN);
  if (rc) return rc;
  const int mt = (g.M + 127) / 128, nt = (g.N + BN - 1) / BN;
  const int nkb = g.K / (fp8 ? 128 : 64);
  int splits = 1;
  const bool plain_f32 = accumulate && g.Cf && !g.Cb && !g.Ct && !g.bias && !g.relu && !g.mask && !g.amaxA;
  /* accumulate: 1 = C is zero already, 2 = zero it here when splitting */
  if (plain_f32) {
    const int sms = ctx().sms > 0 ? ctx().sms : 148;
    while (mt * nt * splits * 2 <= sms && nkb / (splits * 2) >= 8) splits *= 2;
  }
  const int kbps = (nkb + splits - 1) / splits;
  splits = (nkb + kbps - 1) / kbps;
  if (splits > 1 && accumulate == 2) ZCHECK(cudaMemsetAsync(g.Cf, 0, (size_t)g.M * g.N * sizeof(float), s));
  const size_t stage = gemm_stage_bytes(BN);
  if (splits == 1 && (g_gemm_ctas_per_sm == 3 || (g_gemm_ctas_per_sm == 0 && nkb <= kPersistMaxSlices))) {
    /* persistent: a 192 KB ring, one CTA per SM (at least 120 KB of
     * shared memory each, so that two never share an SM's tensor memory) */
    int pst = (int)((192 * 1024) / stage);
    if (pst > kMaxStages) pst = kMaxStages;
    const size_t psmem = std::max<size_t>(1024 + (size_t)pst * stage, 120 * 1024);
    const int sms = ctx().sms > 0 ? ctx().sms : 148;
    const int pgrid = std::min(mt * nt, sms);
#define ZETA_GEMM_PCASE(BNV)                                                                              \
  if (BN == BNV) {                                                                                        \
    auto k = fp8 ? k_gemm_persist<BNV, true> : k_gemm_persist<BNV, false>;                                \
    ZCHECK(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)psmem));              \
    k<<<pgrid, kPersistThreads, psmem, s>>>(ta, tb, g, pst);                                              \
  }
    ZETA_GEMM_PCASE(64)
    ZETA_GEMM_PCASE(128)
    ZETA_GEMM_PCASE(256)
#undef ZETA_GEMM_PCASE
    ZCHECK(cudaGetLastError());
    return ZETA_OK;
  }
  const int ctas = g_gemm_ctas_per_sm == 1 || g_gemm_ctas_per_sm == 2 ? g_gemm_ctas_per_sm : (splits > 1 ? 1 : 2);
  int stages = (int)((ctas == 2 ? 110 * 1024 : 200 * 1024) / stage);
  if (stages > kMaxStages) stages = kMaxStages;
  if (stages > nkb) stages = nkb < 2 ? 2 : nkb;
  const size_t smem = 1024 + (size_t)stages * stage;
  dim3 grid(mt, nt, splits);
#define ZETA_GEMM_CASE(BNV)                                                                              \
  if (BN == BNV) {                                                                                       \
    auto k = fp8 ? k_gemm<BNV, true> : k_gemm<BNV, false>;                                               \
    ZCHECK(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));              \
    k<<<grid, 128, smem, s>>>(ta, tb, g, kbps, stages);                                                  \
  }
  ZETA_GEMM_CASE(64)
  ZETA_GEMM_CASE(128)
  ZETA_GEMM_CASE(256)
#undef ZETA_GEMM_CASE
  ZCHECK(cudaGetLastError());
  return ZETA_OK;
}

}  // namespace zeta

using namespace zeta;

/* Test and tooling entry: C[M x N] (fp32) = A[M x K] . B[N x K]^T with
 * device buffers (bf16, or e4m3 when fp8 != 0).  Returns ZETA_ERR_BUDGET
 * when a tensor-core wait timed out. */
extern "C" int zeta_gemm_configure(int ctas_per_sm) { return gemm_set_ctas_per_sm(ctas_per_sm); }

extern "C" int zeta_gemm_tc(const void *d_A, const void *d_B, float *d_C, int M, int N, int K, int fp8, void *stream) {
  if (!d_A || !d_B || !d_C) return set_error(ZETA_ERR_ARG, "null buffer");
  static uint32_t *d_err = nullptr; /* one error word, kept for the process */
  if (!d_err) ZCHECK(cudaMalloc(&d_err, 4));
  cudaStream_t s = (cudaStream_t)stream;
  ZCHECK(cudaMemsetAsync(d_err, 0, 4, s));
  GemmArgs g{d_A, d_B, M, N, K, nullptr, 0, d_C, nullptr, nullptr, 1.f, d_err, nullptr, nullptr, nullptr};
  int rc = gemm_launch(g, fp8 != 0, s, 2);
  uint32_t err = 0;
  if (rc == ZETA_OK) {
    cudaError_t e = cudaMemcpyAsync(&err, d_err, 4, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) rc = cuda_fail(e, "zeta_gemm_tc");
  }
  if (rc) return rc;
  if (err) return set_error(ZETA_ERR_BUDGET, "gemm: tensor-core wait timed out");
  return ZETA_OK;
}

/* ================================================================== */
/* The network around the GEMMs                                        */
/* ================================================================== */
namespace zeta {
namespace {

constexpr int kIn = 768, kH1 = 512, kH2 = 256, kOut = 128, kEmb = 64;
/* one flat FP32 parameter vector */
constexpr size_t OFF_W1 = 0, OFF_B1 = OFF_W1 + (size_t)kH1 * kIn, OFF_W2 = OFF_B1 + kH1,
                 OFF_B2 = OFF_W2 + (size_t)kH2 * kH1, OFF_W3 = OFF_B2 + kH2, OFF_B3 = OFF_W3 + (size_t)kOut * kH2,
                 OFF_EF = OFF_B3 + kOut, OFF_ET = OFF_EF + (size_t)64 * kEmb, NPARAM = OFF_ET + (size_t)64 * kEmb;
constexpr int kMaxLegal = 218;

/* Input features from the side to move: plane = own/opponent x piece type,
 * square mirrored (sq ^ 56) when black is to move.  Legal moves as
 * (from, to) in the same frame; `target_idx` = index of the target move
 * in that list (-1 when absent or no target given). */
__global__ void k_features(const uint64_t *__restrict__ boards, const uint8_t *__restrict__ stm, const Move *targets,
                           int n, int rows, bf16 *X, bf16 *Xt, uint16_t *moves, uint8_t *nmoves, int16_t *tidx) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= rows) return;
  if (i >= n) { /* padding row: no features, no moves */
    nmoves[i] = 0;
    tidx[i] = -1;
    return;
  }
  const uint64_t *b = boards + 7 * (size_t)i;
  Pos p;
  p.b0 = b[0];
  p.p1 = b[1];
  p.p2 = b[2];
  p.p3 = b[3];
  p.cr = b[4];
  const int s = stm[i] & 1;
  const int flip = s ? 56 : 0;
  u64 occ = p.p1 | p.p2 | p.p3;
  const bf16 one = __float2bfloat16(1.f);
  while (occ) {
    int sq = ctz(occ);
    occ &= occ - 1;
    int pc = piece_at(p, sq);
    int plane = ((pc & 1) != s ? 6 : 0) + (pc >> 1) - 1;
    int f = plane * 64 + (sq ^ flip);
    X[(size_t)i * kIn + f] = one;
    Xt[(size_t)f * rows + i] = one;
  }
  Move list[256];
  int k = gen_legal(p, s, false, list);
  int t = -1;
  const Move target = targets ? (targets[i] & 0x3FFFFFFFu) : 0u;
  for (int j = 0; j < k; j++) {
    Move m = list[j];
    moves[(size_t)i * kMaxLegal + j] = (uint16_t)((m_from(m) ^ flip) | ((m_to(m) ^ flip) << 6));
    if (targets && m == target) t = j;
  }
  nmoves[i] = (uint8_t)k;
  tidx[i] = (int16_t)t;
}

/* Softmax cross-entropy of the legal moves; one warp per position.
 * logit(m) = q_from . Ef[from] + q_to . Et[to].  Writes dQ (and its
 * transpose) scaled by 1/count, accumulates dEf / dEt, the loss and the
 * number of positions whose best-scored move is the target.  With
 * train == 0 it only writes the logits of the moves (scores). */
__global__ void k_head(const float *__restrict__ Q, const float *__restrict__ params, const uint16_t *__restrict__ moves,
                       const uint8_t *__restrict__ nmoves, const int16_t *__restrict__ tidx, int rows, float inv_count,
                       int train, bf16 *dQ, bf16 *dQt, float *grads, float *loss, unsigned *correct, float *scores) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (warp >= rows) return;
  const int i = warp;
  const float *Ef = params + OFF_EF, *Et = params + OFF_ET;
  const float qf0 = Q[(size_t)i * kOut + 2 * lane], qf1 = Q[(size_t)i * kOut + 2 * lane + 1];
  const float qt0 = Q[(size_t)i * kOut + 64 + 2 * lane], qt1 = Q[(size_t)i * kOut + 64 + 2 * lane + 1];
  const int k = nmoves[i];
  const int t = tidx[i];
  /* pass 1: logits (kept in lane j%32, slot j/32) and their maximum */
  float mylog[7];
  float mx = -1e30f;
  int arg = -1;
  for (int j = 0; j < k; j++) {
    const uint16_t mv = moves[(size_t)i * kMaxLegal + j];
    const int f = mv & 63, to = mv >> 6;
    float x = qf0 * Ef[f * 64 + 2 * lane] + qf1 * Ef[f * 64 + 2 * lane + 1] + qt0 * Et[to * 64 + 2 * lane] +
              qt1 * Et[to * 64 + 2 * lane + 1];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xFFFFFFFFu, x, o);
    if ((j & 31) == lane) mylog[j >> 5] = x;
    if (x > mx) {
      mx = x;
      arg = j;
    }
    if (scores) scores[(size_t)i * kMaxLegal + j] = x;
  }
  const int dims[4] = {2 * lane, 2 * lane + 1, 64 + 2 * lane, 64 + 2 * lane + 1};
  if (!train) return;
  if (k == 0 || t < 0) { /* no target: this row adds no gradient */
#pragma unroll
    for (int u = 0; u < 4; u++) {
      dQ[(size_t)i * kOut + dims[u]] = __float2bfloat16(0.f);
      dQt[(size_t)dims[u] * rows + i] = __float2bfloat16(0.f);
    }
    return;
  }
  /* softmax denominator */
  float z = 0.f;
  for (int j = lane; j < k; j += 32) z += __expf(mylog[j >> 5] - mx);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) z += __shfl_xor_sync(0xFFFFFFFFu, z, o);
  const float lt = __shfl_sync(0xFFFFFFFFu, mylog[t >> 5], t & 31);
  if (lane == 0) {
    atomicAdd(loss, (mx + logf(z)) - lt);
    if (arg == t) atomicAdd(correct, 1u);
  }
  /* pass 2: gradients */
  float gf0 = 0.f, gf1 = 0.f, gt0 = 0.f, gt1 = 0.f;
  for (int j = 0; j < k; j++) {
    const float x = __shfl_sync(0xFFFFFFFFu, mylog[j >> 5], j & 31);
    const float dl = (__expf(x - mx) / z - (j == t ? 1.f : 0.f)) * inv_count;
    const uint16_t mv = moves[(size_t)i * kMaxLegal + j];
    const int f = mv & 63, to = mv >> 6;
    gf0 += dl * Ef[f * 64 + 2 * lane];
    gf1 += dl * Ef[f * 64 + 2 * lane + 1];
    gt0 += dl * Et[to * 64 + 2 * lane];
    gt1 += dl * Et[to * 64 + 2 * lane + 1];
    atomicAdd(&grads[OFF_EF + f * 64 + 2 * lane], dl * qf0);
    atomicAdd(&grads[OFF_EF + f * 64 + 2 * lane + 1], dl * qf1);
    atomicAdd(&grads[OFF_ET + to * 64 + 2 * lane], dl * qt0);
    atomicAdd(&grads[OFF_ET + to * 64 + 2 * lane + 1], dl * qt1);
  }
  const float g[4] = {gf0, gf1, gt0, gt1};
#pragma unroll
  for (int u = 0; u < 4; u++) {
    dQ[(size_t)i * kOut + dims[u]] = __float2bfloat16(g[u]);
    dQt[(size_t)dims[u] * rows + i] = __float2bfloat16(g[u]);
  }
}

/* column sums of a rows x cols bf16 matrix into out (bias gradients) */
__global__ void k_colsum(const bf16 *__restrict__ Y, int rows, int cols, float *out) {
  int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= cols) return;
  float s = 0.f;
  for (int r = 0; r < rows; r++) s += __bfloat162float(Y[(size_t)r * cols + c]);
  out[c] = s;
}

/* Adam on the flat parameter vector */
__global__ void k_adam(float *p, const float *g, float *m, float *v, size_t n, float lr, float b1, float b2,
                       float eps, float c1, float c2) {
  size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float gi = g[i];
  float mi = b1 * m[i] + (1.f - b1) * gi, vi = b2 * v[i] + (1.f - b2) * gi * gi;
  m[i] = mi;
  v[i] = vi;
  p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
}

/* BF16 copies of a rows x cols FP32 weight: as is, and transposed */
__global__ void k_to_bf16(const float *__restrict__ W, int rows, int cols, bf16 *Wb, bf16 *Wt) {
  size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (size_t)rows * cols) return;
  int r = (int)(i / cols), c = (int)(i % cols);
  bf16 x = __float2bfloat16(W[i]);
  if (Wb) Wb[i] = x;
  if (Wt) Wt[(size_t)c * rows + r] = x;
}

/* FP8 E4M3 copy with a per-tensor scale: q = x / scale, scale = max|x|/448 */
__global__ void k_absmax(const float *__restrict__ x, size_t n, unsigned *out_bits) {
  size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  float a = i < n ? fabsf(x[i]) : 0.f;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) a = fmaxf(a, __shfl_xor_sync(0xFFFFFFFFu, a, o));
  if ((threadIdx.x & 31) == 0) atomicMax(out_bits, __float_as_uint(a)); /* non-negative floats order as ints */
}
__global__ void k_absmax_bf16(const bf16 *__restrict__ x, size_t n, unsigned *out_bits) {
  size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  float a = i < n ? fabsf(__bfloat162float(x[i])) : 0.f;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) a = fmaxf(a, __shfl_xor_sync(0xFFFFFFFFu, a, o));
  if ((threadIdx.x & 31) == 0) atomicMax(out_bits, __float_as_uint(a));
}
__global__ void k_quant_fp8(const float *__restrict__ xf, const bf16 *__restrict__ xb, size_t n,
                            const unsigned *absmax_bits, __nv_fp8_e4m3 *q) {
  size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float am = __uint_as_float(*absmax_bits);
  float inv = am > 0.f ? 448.f / am : 1.f;
  float x = xf ? xf[i] : __bfloat162float(xb[i]);
  q[i] = __nv_fp8_e4m3(x * inv);
}

/* ---------------- state ---------------- */
struct MlpState {
  float *params = nullptr, *grads = nullptr, *m = nullptr, *v = nullptr;
  bf16 *W1b = nullptr, *W2b = nullptr, *W3b = nullptr, *W2t = nullptr, *W3t = nullptr;
  __nv_fp8_e4m3 *W1q = nullptr, *W2q = nullptr, *W3q = nullptr;
  unsigned *amax = nullptr; /* [0..2] weights, [3..5] activations (float bits) */
  int cap = 0;              /* activation rows */
  bf16 *X = nullptr, *Xt = nullptr, *H1 = nullptr, *H1t = nullptr, *H2 = nullptr, *H2t = nullptr;
  bf16 *dQ = nullptr, *dQt = nullptr, *dH2 = nullptr, *dH2t = nullptr, *dH1 = nullptr, *dH1t = nullptr;
  __nv_fp8_e4m3 *Xq = nullptr, *H1q = nullptr, *H2q = nullptr;
  float *Q = nullptr, *scores = nullptr;
  uint16_t *moves = nullptr;
  uint8_t *nmoves = nullptr;
  int16_t *tidx = nullptr;
  float *loss = nullptr;
  unsigned *correct = nullptr;
  uint32_t *err = nullptr;
  uint64_t *d_boards = nullptr;
  uint8_t *d_stm = nullptr;
  Move *d_targets = nullptr;
  int data_cap = 0;
  int step = 0;
};

MlpState *state() { return (MlpState *)ctx().mlp; }

unsigned long long g_rng;
float urand() { /* splitmix64 -> [0,1) */
  unsigned long long z = (g_rng += 0x9E3779B97F4A7C15ULL);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  z ^= z >> 31;
  return (float)((z >> 11) * (1.0 / 9007199254740992.0));
}

template <typename T>
int dalloc(T *&p, size_t n) {
  ZCHECK(cudaMalloc(&p, n * sizeof(T)));
  return ZETA_OK;
}

int ensure_rows(MlpState &S, int rows) {
  if (rows <= S.cap) return ZETA_OK;
  void *bufs[] = {S.X, S.Xt, S.H1, S.H1t, S.H2, S.H2t, S.dQ, S.dQt, S.dH2, S.dH2t, S.dH1, S.dH1t,
                  S.Xq, S.H1q, S.H2q, S.Q, S.scores, S.moves, S.nmoves, S.tidx};
  for (void *b : bufs) cudaFree(b);
  const size_t R = (size_t)rows;
  int rc = 0;
  rc |= dalloc(S.X, R * kIn) | dalloc(S.Xt, R * kIn) | dalloc(S.H1, R * kH1) | dalloc(S.H1t, R * kH1);
  rc |= dalloc(S.H2, R * kH2) | dalloc(S.H2t, R * kH2) | dalloc(S.dQ, R * kOut) | dalloc(S.dQt, R * kOut);
  rc |= dalloc(S.dH2, R * kH2) | dalloc(S.dH2t, R * kH2) | dalloc(S.dH1, R * kH1) | dalloc(S.dH1t, R * kH1);
  rc |= dalloc(S.Xq, R * kIn) | dalloc(S.H1q, R * kH1) | dalloc(S.H2q, R * kH2) | dalloc(S.Q, R * kOut);
  rc |= dalloc(S.scores, R * kMaxLegal) | dalloc(S.moves, R * kMaxLegal) | dalloc(S.nmoves, R) | dalloc(S.tidx, R);
  if (rc) return ZETA_ERR_CUDA;
  S.cap = rows;
  return ZETA_OK;
}

/* BF16 and FP8 copies of the weights after every update */
int refresh_weights(MlpState &S, cudaStream_t s) {
  auto grid = [](size_t n) { return (unsigned)((n + 255) / 256); };
  k_to_bf16<<<grid((size_t)kH1 * kIn), 256, 0, s>>>(S.params + OFF_W1, kH1, kIn, S.W1b, nullptr);
  k_to_bf16<<<grid((size_t)kH2 * kH1), 256, 0, s>>>(S.params + OFF_W2, kH2, kH1, S.W2b, S.W2t);
  k_to_bf16<<<grid((size_t)kOut * kH2), 256, 0, s>>>(S.params + OFF_W3, kOut, kH2, S.W3b, S.W3t);
  ZCHECK(cudaMemsetAsync(S.amax, 0, 3 * sizeof(unsigned), s));
  const size_t off[3] = {OFF_W1, OFF_W2, OFF_W3}, num[3] = {(size_t)kH1 * kIn, (size_t)kH2 * kH1, (size_t)kOut * kH2};
  __nv_fp8_e4m3 *q[3] = {S.W1q, S.W2q, S.W3q};
  for (int i = 0; i < 3; i++) {
    k_absmax<<<grid(num[i]), 256, 0, s>>>(S.params + off[i], num[i], S.amax + i);
    k_quant_fp8<<<grid(num[i]), 256, 0, s>>>(S.params + off[i], nullptr, num[i], S.amax + i, q[i]);
  }
  ZCHECK(cudaGetLastError());
  return ZETA_OK;
}

int mlp_create(unsigned long long seed) {
  Context &c = ctx();
  if (!c.mlp) c.mlp = new MlpState();
  MlpState &S = *state();
  if (!S.params) {
    int rc = dalloc(S.params, NPARAM) | dalloc(S.grads, NPARAM) | dalloc(S.m, NPARAM) | dalloc(S.v, NPARAM);
    rc |= dalloc(S.W1b, (size_t)kH1 * kIn) | dalloc(S.W2b, (size_t)kH2 * kH1) | dalloc(S.W3b, (size_t)kOut * kH2);
    rc |= dalloc(S.W2t, (size_t)kH2 * kH1) | dalloc(S.W3t, (size_t)kOut * kH2);
    rc |= dalloc(S.W1q, (size_t)kH1 * kIn) | dalloc(S.W2q, (size_t)kH2 * kH1) | dalloc(S.W3q, (size_t)kOut * kH2);
    rc |= dalloc(S.amax, 8) | dalloc(S.loss, 1) | dalloc(S.correct, 1) | dalloc(S.err, 1);
    if (rc) return ZETA_ERR_CUDA;
  }
  /* He-uniform weights, zero biases, small embeddings */
  std::vector<float> h(NPARAM, 0.f);
  g_rng = seed;
  auto fill = [&](size_t off, size_t n, float lim) {
    for (size_t i = 0; i < n; i++) h[off + i] = (2.f * urand() - 1.f) * lim;
  };
  fill(OFF_W1, (size_t)kH1 * kIn, sqrtf(6.f / 32.f)); /* about 32 active inputs */
  fill(OFF_W2, (size_t)kH2 * kH1, sqrtf(6.f / kH1));
  fill(OFF_W3, (size_t)kOut * kH2, sqrtf(3.f / kH2));
  fill(OFF_EF, (size_t)64 * kEmb, 0.5f);
  fill(OFF_ET, (size_t)64 * kEmb, 0.5f);
  ZCHECK(cudaMemcpy(S.params, h.data(), NPARAM * sizeof(float), cudaMemcpyHostToDevice));
  ZCHECK(cudaMemset(S.m, 0, NPARAM * sizeof(float)));
  ZCHECK(cudaMemset(S.v, 0, NPARAM * sizeof(float)));
  S.step = 0;
  int rc = refresh_weights(S, c.stream);
  if (rc) return rc;
  ZCHECK(cudaStreamSynchronize(c.stream));
  return ZETA_OK;
}

GemmArgs gemm(const void *A, const void *B, int M, int N, int K, uint32_t *err) {
  GemmArgs g{A, B, M, N, K, nullptr, 0, nullptr, nullptr, nullptr, 1.f, err, nullptr, nullptr, nullptr};
  return g;
}

/* features, move lists and the forward pass of `rows` positions
 * (rows a multiple of 128; n real ones) */
int forward(MlpState &S, const uint64_t *d_boards, const uint8_t *d_stm, const Move *d_targets, int n, int rows,
            bool fp8, cudaStream_t s) {
  int rc;
  ZCHECK(cudaMemsetAsync(S.X, 0, (size_t)rows * kIn * sizeof(bf16), s));
  ZCHECK(cudaMemsetAsync(S.Xt, 0, (size_t)rows * kIn * sizeof(bf16), s));
  k_features<<<(rows + 127) / 128, 128, 0, s>>>(d_boards, d_stm, d_targets, n, rows, S.X, S.Xt, S.moves, S.nmoves,
                                                S.tidx);
  ZCHECK(cudaGetLastError());
  const float *P = S.params;
  if (!fp8) {
    GemmArgs g1 = gemm(S.X, S.W1b, rows, kH1, kIn, S.err);
    g1.bias = P + OFF_B1, g1.relu = 1, g1.Cb = S.H1, g1.Ct = S.H1t;
    if ((rc = gemm_launch(g1, false, s))) return rc;
    GemmArgs g2 = gemm(S.H1, S.W2b, rows, kH2, kH1, S.err);
    g2.bias = P + OFF_B2, g2.relu = 1, g2.Cb = S.H2, g2.Ct = S.H2t;
    if ((rc = gemm_launch(g2, false, s))) return rc;
    GemmArgs g3 = gemm(S.H2, S.W3b, rows, kOut, kH2, S.err);
    g3.bias = P + OFF_B3, g3.Cf = S.Q;
    return gemm_launch(g3, false, s);
  }
  /* FP8 E4M3 inference: per-tensor scales of the activations, measured */
  auto grid = [](size_t n) { return (unsigned)((n + 255) / 256); };
  ZCHECK(cudaMemsetAsync(S.amax + 3, 0, 3 * sizeof(unsigned), s));
  size_t nx = (size_t)rows * kIn;
  k_absmax_bf16<<<grid(nx), 256, 0, s>>>(S.X, nx, S.amax + 3);
  k_quant_fp8<<<grid(nx), 256, 0, s>>>(nullptr, S.X, nx, S.amax + 3, S.Xq);
  GemmArgs g1 = gemm(S.Xq, S.W1q, rows, kH1, kIn, S.err);
  g1.bias = P + OFF_B1, g1.relu = 1, g1.Cb = S.H1, g1.amaxA = S.amax + 3, g1.amaxB = S.amax + 0;
  if ((rc = gemm_launch(g1, true, s))) return rc;
  size_t nh1 = (size_t)rows * kH1;
  k_absmax_bf16<<<grid(nh1), 256, 0, s>>>(S.H1, nh1, S.amax + 4);
  k_quant_fp8<<<grid(nh1), 256, 0, s>>>(nullptr, S.H1, nh1, S.amax + 4, S.H1q);
  GemmArgs g2 = gemm(S.H1q, S.W2q, rows, kH2, kH1, S.err);
  g2.bias = P + OFF_B2, g2.relu = 1, g2.Cb = S.H2, g2.amaxA = S.amax + 4, g2.amaxB = S.amax + 1;
  if ((rc = gemm_launch(g2, true, s))) return rc;
  size_t nh2 = (size_t)rows * kH2;
  k_absmax_bf16<<<grid(nh2), 256, 0, s>>>(S.H2, nh2, S.amax + 5);
  k_quant_fp8<<<grid(nh2), 256, 0, s>>>(nullptr, S.H2, nh2, S.amax + 5, S.H2q);
  GemmArgs g3 = gemm(S.H2q, S.W3q, rows, kOut, kH2, S.err);
  g3.bias = P + OFF_B3, g3.Cf = S.Q, g3.amaxA = S.amax + 5, g3.amaxB = S.amax + 2;
  return gemm_launch(g3, true, s);
}

/* loss head and the backward pass into S.grads (mean over n positions) */
int backward(MlpState &S, int n, int rows, cudaStream_t s) {
  int rc;
  ZCHECK(cudaMemsetAsync(S.grads, 0, NPARAM * sizeof(float), s));
  k_head<<<(rows * 32 + 127) / 128, 128, 0, s>>>(S.Q, S.params, S.moves, S.nmoves, S.tidx, rows, 1.f / (float)n, 1,
                                                 S.dQ, S.dQt, S.grads, S.loss, S.correct, nullptr);
  ZCHECK(cudaGetLastError());
  float *G = S.grads;
  GemmArgs a = gemm(S.dQ, S.W3t, rows, kH2, kOut, S.err); /* dH2 = dQ W3 . relu'(H2) */
  a.mask = S.H2, a.Cb = S.dH2, a.Ct = S.dH2t;
  if ((rc = gemm_launch(a, false, s))) return rc;
  GemmArgs b = gemm(S.dQt, S.H2t, kOut, kH2, rows, S.err); /* dW3 = dQ^T H2 */
  b.Cf = G + OFF_W3;
  if ((rc = gemm_launch(b, false, s, 1))) return rc; /* into the zeroed gradient */
  GemmArgs c = gemm(S.dH2, S.W2t, rows, kH1, kH2, S.err); /* dH1 = dH2 W2 . relu'(H1) */
  c.mask = S.H1, c.Cb = S.dH1, c.Ct = S.dH1t;
  if ((rc = gemm_launch(c, false, s))) return rc;
  GemmArgs d = gemm(S.dH2t, S.H1t, kH2, kH1, rows, S.err); /* dW2 = dH2^T H1 */
  d.Cf = G + OFF_W2;
  if ((rc = gemm_launch(d, false, s, 1))) return rc; /* into the zeroed gradient */
  GemmArgs e = gemm(S.dH1t, S.Xt, kH1, kIn, rows, S.err); /* dW1 = dH1^T X */
  e.Cf = G + OFF_W1;
  if ((rc = gemm_launch(e, false, s, 1))) return rc; /* into the zeroed gradient */
  k_colsum<<<(kOut + 127) / 128, 128, 0, s>>>(S.dQ, rows, kOut, G + OFF_B3);
  k_colsum<<<(kH2 + 127) / 128, 128, 0, s>>>(S.dH2, rows, kH2, G + OFF_B2);
  k_colsum<<<(kH1 + 127) / 128, 128, 0, s>>>(S.dH1, rows, kH1, G + OFF_B1);
  ZCHECK(cudaGetLastError());
  return ZETA_OK;
}

int load_data(MlpState &S, const uint64_t *boards, const uint8_t *stm, const uint32_t *targets, int n,
              cudaStream_t s) {
  if (n > S.data_cap) {
    cudaFree(S.d_boards);
    cudaFree(S.d_stm);
    cudaFree(S.d_targets);
    S.data_cap = 0;
    int rc = dalloc(S.d_boards, (size_t)n * 7) | dalloc(S.d_stm, (size_t)n) | dalloc(S.d_targets, (size_t)n);
    if (rc) return ZETA_ERR_CUDA;
    S.data_cap = n;
  }
  ZCHECK(cudaMemcpyAsync(S.d_boards, boards, (size_t)n * 56, cudaMemcpyHostToDevice, s));
  ZCHECK(cudaMemcpyAsync(S.d_stm, stm, (size_t)n, cudaMemcpyHostToDevice, s));
  if (targets) ZCHECK(cudaMemcpyAsync(S.d_targets, targets, (size_t)n * 4, cudaMemcpyHostToDevice, s));
  return ZETA_OK;
}

/* search requests -> board rows for the feature kernel */
__global__ void k_req_to_boards(const OrderRequest *__restrict__ req, int n, uint64_t *boards, uint8_t *stm) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const OrderRequest q = req[i];
  uint64_t *b = boards + 7 * (size_t)i;
  for (int k = 0; k < 5; k++) b[k] = q.b[k];
  b[5] = q.key;
  b[6] = 0;
  stm[i] = (uint8_t)q.stm;
}

/* the 12 highest-scored moves of each row into the ordering cache, as
 * real-board (from | to << 6) */
__global__ void k_topk_cache(const OrderRequest *__restrict__ req, int n, const float *__restrict__ scores,
                             const uint16_t *__restrict__ moves, const uint8_t *__restrict__ nmoves, OrderEntry *cache,
                             unsigned long long mask) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int k = nmoves[i];
  const int flip = req[i].stm ? 56 : 0;
  float bs[kOrderTop];
  int bi[kOrderTop];
#pragma unroll
  for (int r = 0; r < kOrderTop; r++) {
    bs[r] = -1e30f;
    bi[r] = -1;
  }
  for (int j = 0; j < k; j++) {
    float x = scores[(size_t)i * kMaxLegal + j];
    if (x <= bs[kOrderTop - 1]) continue;
    int r = kOrderTop - 1;
    while (r > 0 && bs[r - 1] < x) {
      bs[r] = bs[r - 1];
      bi[r] = bi[r - 1];
      r--;
    }
    bs[r] = x;
    bi[r] = j;
  }
  OrderEntry e;
  e.key = req[i].key;
#pragma unroll
  for (int r = 0; r < kOrderTop; r++) {
    if (bi[r] < 0) {
      e.mv[r] = 0xFFFF;
    } else {
      const uint16_t mv = moves[(size_t)i * kMaxLegal + bi[r]];
      e.mv[r] = (uint16_t)(((mv & 63) ^ flip) | ((((mv >> 6) & 63) ^ flip) << 6));
    }
  }
  cache[e.key & mask] = e;
}

int ensure_data(MlpState &S, int n) {
  if (n <= S.data_cap) return ZETA_OK;
  cudaFree(S.d_boards);
  cudaFree(S.d_stm);
  cudaFree(S.d_targets);
  S.data_cap = 0;
  int rc = dalloc(S.d_boards, (size_t)n * 7) | dalloc(S.d_stm, (size_t)n) | dalloc(S.d_targets, (size_t)n);
  if (rc) return ZETA_ERR_CUDA;
  S.data_cap = n;
  return ZETA_OK;
}

int check_err(MlpState &S, cudaStream_t s) {
  uint32_t e = 0;
  ZCHECK(cudaMemcpyAsync(&e, S.err, 4, cudaMemcpyDeviceToHost, s));
  ZCHECK(cudaStreamSynchronize(s));
  if (e) return set_error(ZETA_ERR_BUDGET, "mlp: a tensor-core wait timed out");
  return ZETA_OK;
}

}  // namespace

bool mlp_ready_for_search() { return ctx().mlp && state()->params; }

int mlp_fill_order_cache(const OrderRequest *req, uint32_t nreq, OrderEntry *cache, uint64_t mask, int fp8,
                         cudaStream_t s) {
  MlpState &S = *state();
  const int chunk = 16384;
  int rc;
  if ((rc = ensure_rows(S, chunk)) || (rc = ensure_data(S, chunk))) return rc;
  ZCHECK(cudaMemsetAsync(S.err, 0, 4, s));
  for (uint32_t off = 0; off < nreq; off += chunk) {
    const int cnt = (int)(nreq - off < (uint32_t)chunk ? nreq - off : (uint32_t)chunk);
    const int rows = (cnt + 127) / 128 * 128;
    k_req_to_boards<<<(cnt + 127) / 128, 128, 0, s>>>(req + off, cnt, S.d_boards, S.d_stm);
    ZCHECK(cudaGetLastError());
    if ((rc = forward(S, S.d_boards, S.d_stm, nullptr, cnt, rows, fp8 != 0, s))) return rc;
    k_head<<<(rows * 32 + 127) / 128, 128, 0, s>>>(S.Q, S.params, S.moves, S.nmoves, S.tidx, rows, 1.f, 0, nullptr,
                                                   nullptr, nullptr, nullptr, nullptr, S.scores);
    k_topk_cache<<<(cnt + 127) / 128, 128, 0, s>>>(req + off, cnt, S.scores, S.moves, S.nmoves, cache, mask);
    ZCHECK(cudaGetLastError());
  }
  return check_err(S, s);
}

void mlp_free() {
  Context &c = ctx();
  MlpState *S = (MlpState *)c.mlp;
  if (!S) return;
  void *bufs[] = {S->params, S->grads, S->m, S->v, S->W1b, S->W2b, S->W3b, S->W2t, S->W3t, S->W1q, S->W2q,
                  S->W3q, S->amax, S->X, S->Xt, S->H1, S->H1t, S->H2, S->H2t, S->dQ, S->dQt, S->dH2, S->dH2t,
                  S->dH1, S->dH1t, S->Xq, S->H1q, S->H2q, S->Q, S->scores, S->moves, S->nmoves, S->tidx,
                  S->loss, S->correct, S->err, S->d_boards, S->d_stm, S->d_targets};
  for (void *b : bufs) cudaFree(b);
  delete S;
  c.mlp = nullptr;
}

}  // namespace zeta

static int mlp_ready() {
  if (!zeta::ctx().ready) return set_error(ZETA_ERR_STATE, "zeta_init has not been called");
  if (!zeta::ctx().mlp || !((zeta::MlpState *)zeta::ctx().mlp)->params)
    return set_error(ZETA_ERR_STATE, "zeta_mlp_init has not been called");
  return ZETA_OK;
}

extern "C" {

int zeta_mlp_init(uint64_t seed) {
  if (!ctx().ready) return set_error(ZETA_ERR_STATE, "zeta_init has not been called");
  return mlp_create(seed);
}

int zeta_mlp_param_count(void) { return (int)NPARAM; }

int zeta_mlp_get_params(float *out) {
  int rc = mlp_ready();
  if (rc) return rc;
  ZCHECK(cudaMemcpy(out, state()->params, NPARAM * sizeof(float), cudaMemcpyDeviceToHost));
  return ZETA_OK;
}

int zeta_mlp_set_params(const float *in) {
  int rc = mlp_ready();
  if (rc) return rc;
  MlpState &S = *state();
  ZCHECK(cudaMemcpy(S.params, in, NPARAM * sizeof(float), cudaMemcpyHostToDevice));
  rc = refresh_weights(S, ctx().stream);
  if (rc) return rc;
  ZCHECK(cudaStreamSynchronize(ctx().stream));
  return ZETA_OK;
}

/* One batch: forward, loss and gradients (no update).  grads: NPARAM
 * floats in the flat layout of zeta_mlp_get_params; loss: mean. */
int zeta_mlp_grads(const uint64_t *boards, const uint8_t *stm, const uint32_t *targets, int n, float *grads,
                   float *loss) {
  int rc = mlp_ready();
  if (rc) return rc;
  if (n <= 0) return set_error(ZETA_ERR_ARG, "empty batch");
  MlpState &S = *state();
  cudaStream_t s = ctx().stream;
  const int rows = (n + 127) / 128 * 128;
  if ((rc = ensure_rows(S, rows)) || (rc = load_data(S, boards, stm, targets, n, s))) return rc;
  ZCHECK(cudaMemsetAsync(S.err, 0, 4, s));
  ZCHECK(cudaMemsetAsync(S.loss, 0, 4, s));
  ZCHECK(cudaMemsetAsync(S.correct, 0, 4, s));
  if ((rc = forward(S, S.d_boards, S.d_stm, S.d_targets, n, rows, false, s))) return rc;
  if ((rc = backward(S, n, rows, s))) return rc;
  if ((rc = check_err(S, s))) return rc;
  if (grads) ZCHECK(cudaMemcpy(grads, S.grads, NPARAM * sizeof(float), cudaMemcpyDeviceToHost));
  float l = 0;
  ZCHECK(cudaMemcpy(&l, S.loss, 4, cudaMemcpyDeviceToHost));
  if (loss) *loss = l / (float)n;
  return ZETA_OK;
}

/* Adam training over (boards, stm, best move) examples, `epochs` passes in
 * order, batches of `batch` (a multiple of 128).  Per epoch: mean loss
 * and the share of examples whose highest-scored legal move is the
 * target (the model's state before each update). */
int zeta_mlp_train(const uint64_t *boards, const uint8_t *stm, const uint32_t *targets, int n, int epochs, int batch,
                   float lr, float *loss_per_epoch, float *acc_per_epoch) {
  int rc = mlp_ready();
  if (rc) return rc;
  if (n <= 0 || epochs <= 0 || batch <= 0 || batch % 128) return set_error(ZETA_ERR_ARG, "bad training arguments");
  MlpState &S = *state();
  cudaStream_t s = ctx().stream;
  if ((rc = ensure_rows(S, batch)) || (rc = load_data(S, boards, stm, targets, n, s))) return rc;
  ZCHECK(cudaMemsetAsync(S.err, 0, 4, s));
  const float b1 = 0.9f, b2 = 0.999f;
  for (int ep = 0; ep < epochs; ep++) {
    ZCHECK(cudaMemsetAsync(S.loss, 0, 4, s));
    ZCHECK(cudaMemsetAsync(S.correct, 0, 4, s));
    for (int off = 0; off < n; off += batch) {
      const int cnt = n - off < batch ? n - off : batch;
      const int rows = (cnt + 127) / 128 * 128;
      if ((rc = forward(S, S.d_boards + 7 * (size_t)off, S.d_stm + off, S.d_targets + off, cnt, rows, false, s)))
        return rc;
      if ((rc = backward(S, cnt, rows, s))) return rc;
      S.step++;
      const float c1 = 1.f - powf(b1, (float)S.step), c2 = 1.f - powf(b2, (float)S.step);
      k_adam<<<(unsigned)((NPARAM + 255) / 256), 256, 0, s>>>(S.params, S.grads, S.m, S.v, NPARAM, lr, b1, b2, 1e-8f,
                                                             c1, c2);
      ZCHECK(cudaGetLastError());
      if ((rc = refresh_weights(S, s))) return rc;
    }
    float l = 0;
    unsigned corr = 0;
    ZCHECK(cudaMemcpyAsync(&l, S.loss, 4, cudaMemcpyDeviceToHost, s));
    ZCHECK(cudaMemcpyAsync(&corr, S.correct, 4, cudaMemcpyDeviceToHost, s));
    if ((rc = check_err(S, s))) return rc;
    if (loss_per_epoch) loss_per_epoch[ep] = l / (float)n;
    if (acc_per_epoch) acc_per_epoch[ep] = (float)corr / (float)n;
  }
  return ZETA_OK;
}

/* Scores of every legal move of n positions (BF16, or FP8 E4M3 when fp8 !=
 * 0): scores n x 218 floats in the order of the engine's move generator,
 * nmoves n counts; the engine orders by them.  best (optional): index of
 * the highest score. */
int zeta_mlp_scores(const uint64_t *boards, const uint8_t *stm, int n, int fp8, float *scores, uint8_t *nmoves,
                    int32_t *best) {
  int rc = mlp_ready();
  if (rc) return rc;
  if (n <= 0) return set_error(ZETA_ERR_ARG, "empty batch");
  MlpState &S = *state();
  cudaStream_t s = ctx().stream;
  const int rows = (n + 127) / 128 * 128;
  if ((rc = ensure_rows(S, rows)) || (rc = load_data(S, boards, stm, nullptr, n, s))) return rc;
  ZCHECK(cudaMemsetAsync(S.err, 0, 4, s));
  if ((rc = forward(S, S.d_boards, S.d_stm, nullptr, n, rows, fp8 != 0, s))) return rc;
  k_head<<<(rows * 32 + 127) / 128, 128, 0, s>>>(S.Q, S.params, S.moves, S.nmoves, S.tidx, rows, 1.f, 0, nullptr,
                                                 nullptr, nullptr, nullptr, nullptr, S.scores);
  ZCHECK(cudaGetLastError());
  if ((rc = check_err(S, s))) return rc;
  std::vector<float> sc((size_t)n * kMaxLegal);
  std::vector<uint8_t> nm(n);
  ZCHECK(cudaMemcpy(sc.data(), S.scores, sc.size() * 4, cudaMemcpyDeviceToHost));
  ZCHECK(cudaMemcpy(nm.data(), S.nmoves, n, cudaMemcpyDeviceToHost));
  if (scores) memcpy(scores, sc.data(), sc.size() * 4);
  if (nmoves) memcpy(nmoves, nm.data(), n);
  if (best)
    for (int i = 0; i < n; i++) {
      int b = -1;
      float bv = -1e30f;
      for (int j = 0; j < nm[i]; j++)
        if (sc[(size_t)i * kMaxLegal + j] > bv) bv = sc[(size_t)i * kMaxLegal + j], b = j;
      best[i] = b;
    }
  return ZETA_OK;
}

}  // extern "C"
