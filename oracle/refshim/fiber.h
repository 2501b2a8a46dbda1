/*
 * fiber.h -- 64-lane work-group emulator for the reference kernels
 * (TEST INFRASTRUCTURE ONLY).  Portable C/C++: ucontext creates each
 * fiber's stack once; switches are _setjmp/_longjmp, which avoid the
 * signal-mask system call of swapcontext.  No inline assembly, so the same
 * source builds on x86-64 and aarch64.
 */
#ifndef REFSHIM_FIBER_H
#define REFSHIM_FIBER_H

namespace refshim {

/* Run body(arg) as `lanes` fibers on the calling thread until every fiber
 * returns.  The body must execute the same number of barriers per lane
 * (true of both reference kernels). */
void run_workgroup(void (*body)(void *), void *arg, int lanes);

/* Lane id of the running fiber. */
int fiber_lane();

/* Work-group barrier: switch to the next lane. */
void fiber_yield();

/* global ids 0/1 and sizes 0/1 reported to the kernel running on this thread */
void set_work_item(unsigned long id0, unsigned long id1, unsigned long size0, unsigned long size1);

}  // namespace refshim

#endif
