/*
 * peak.cu -- integer-ALU throughput of the GPU, measured.
 *
 * The perft and search kernels are bound by 32-bit logic, shift and add
 * instructions (every u64 bitboard operation is two of them).  No
 * datasheet figure is used: this kernel issues only lop3.b32 and
 * shf.l.wrap.b32 (the instructions the bitboard code compiles to) in 8
 * independent chains per thread on every SM and reports operations per
 * second, one operation per 32-bit instruction per thread.
 */
#include "context.cuh"

namespace zeta {

namespace {
constexpr int kChains = 8;
constexpr int kIters = 4096;

__global__ void __launch_bounds__(256) k_int_peak(uint32_t seed, uint32_t *out) {
  uint32_t a[kChains], b[kChains];
#pragma unroll
  for (int c = 0; c < kChains; c++) {
    a[c] = seed ^ (threadIdx.x * 0x9E3779B9u + c);
    b[c] = seed + blockIdx.x * 977u + c * 131u;
  }
  for (int i = 0; i < kIters; i++) {
#pragma unroll
    for (int c = 0; c < kChains; c++) {
      asm volatile("lop3.b32 %0, %0, %1, %2, 0x96;" : "+r"(a[c]) : "r"(b[c]), "r"(seed));
      asm volatile("shf.l.wrap.b32 %0, %0, %1, 7;" : "+r"(b[c]) : "r"(a[c]));
    }
  }
  uint32_t x = 0;
#pragma unroll
  for (int c = 0; c < kChains; c++) x ^= a[c] ^ b[c];
  if (x == 0x12345678u) out[0] = x; /* keeps the chains live */
}
}  // namespace

int int_peak(double *tops) {
  Context &c = ctx();
  uint32_t *d_out = nullptr;
  ZCHECK(cudaMalloc(&d_out, 4));
  int bps = 0;
  ZCHECK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, k_int_peak, 256, 0));
  int blocks = c.sms * (bps > 0 ? bps : 1);
  for (int w = 0; w < 2; w++) k_int_peak<<<blocks, 256, 0, c.stream>>>(1u + w, d_out);
  ZCHECK(cudaGetLastError());
  ZCHECK(cudaEventRecord(c.ev[0], c.stream));
  const int reps = 5;
  for (int r = 0; r < reps; r++) k_int_peak<<<blocks, 256, 0, c.stream>>>(7u + r, d_out);
  ZCHECK(cudaEventRecord(c.ev[1], c.stream));
  ZCHECK(cudaEventSynchronize(c.ev[1]));
  float ms = 0;
  ZCHECK(cudaEventElapsedTime(&ms, c.ev[0], c.ev[1]));
  cudaFree(d_out);
  double ops = (double)reps * blocks * 256.0 * kIters * kChains * 2.0;
  *tops = ops / (ms * 1e-3) / 1e12;
  return ZETA_OK;
}

}  // namespace zeta
