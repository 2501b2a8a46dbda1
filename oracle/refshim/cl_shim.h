/*
 * cl_shim.h -- maps the OpenCL C dialect used by the reference kernels
 * (src/zetaperft.cl, src/zeta.cl) onto C++ so that the unmodified kernel
 * sources compile as host code.  TEST INFRASTRUCTURE ONLY (oracle).
 *
 * One work-group of 64 work-items becomes 64 fibers on one OS thread
 * (fiber.h); barrier() switches to the next fiber, so a barrier phase runs
 * lanes 0..63 in order.  __local variables are thread_local statics, shared
 * by the fibers of the work-group that the thread is running.
 * __OPENCL_VERSION__ stays undefined, which selects the kernels' SWAR
 * popcount and their serial (OLDSCHOOL) reductions: both deterministic.
 */
#ifndef REFSHIM_CL_SHIM_H
#define REFSHIM_CL_SHIM_H

#include "fiber.h"

/* no system headers: this file is preprocessed on one machine and may be
 * compiled on another (x86-64 here, aarch64 on the GPU host) */
typedef __SIZE_TYPE__ size_t;

typedef unsigned long ulong;
typedef unsigned int uint;
typedef unsigned char uchar;

#define __kernel
#define __global
#define __private
#define __constant static const
#define __local static thread_local

#define CLK_LOCAL_MEM_FENCE 1
#define CLK_GLOBAL_MEM_FENCE 2

namespace refshim {
/* work-item ids of the running fiber */
struct WorkItem {
  size_t global_id[3];
  size_t global_size[3];
};
extern thread_local WorkItem g_item;
}  // namespace refshim

static inline void barrier(int) { refshim::fiber_yield(); }
static inline size_t get_local_id(int d) { return d == 2 ? (size_t)refshim::fiber_lane() : 0; }
static inline size_t get_global_id(int d) {
  return d == 2 ? (size_t)refshim::fiber_lane() : refshim::g_item.global_id[d];
}
static inline size_t get_global_size(int d) { return d == 2 ? 64 : refshim::g_item.global_size[d]; }

/* OpenCL atomics on global memory: real atomics, so work-groups running on
 * several OS threads (ABDADA workers) share the tables correctly. */
template <class T, class A, class B>
static inline T atom_cmpxchg(T *p, A cmp, B val) {
  T expected = (T)cmp;
  __atomic_compare_exchange_n(p, &expected, (T)val, false, __ATOMIC_SEQ_CST, __ATOMIC_SEQ_CST);
  return expected;
}
template <class T, class A>
static inline T atom_xchg(T *p, A val) {
  return __atomic_exchange_n(p, (T)val, __ATOMIC_SEQ_CST);
}

#endif
