/*
 * fiber.cc -- work-group emulator (see fiber.h).  TEST INFRASTRUCTURE ONLY.
 */
#include "fiber.h"

#include <setjmp.h>
#include <stdio.h>
#include <stdlib.h>
#include <ucontext.h>

#include "cl_shim.h"

namespace refshim {

thread_local WorkItem g_item = {{0, 0, 0}, {1, 1, 64}};

namespace {
constexpr int kMaxLanes = 64;
constexpr size_t kStack = 256 * 1024;

struct Lane {
  jmp_buf ctx;
  ucontext_t boot;
  char *stack;
  bool done;
};

struct Group {
  Lane lane[kMaxLanes];
  int nlanes;
  int cur;
  jmp_buf sched;
  ucontext_t sched_uc;
  void (*body)(void *);
  void *arg;
};

thread_local Group *g_group = nullptr;

void trampoline() {
  Group *g = g_group;
  int id = g->cur;
  /* park: record this lane's entry point and return to the scheduler */
  if (_setjmp(g->lane[id].ctx) == 0) _longjmp(g->sched, 1);
  g = g_group;
  g->body(g->arg);
  g->lane[g->cur].done = true;
  _longjmp(g->sched, 1);
}
}  // namespace

void set_work_item(unsigned long id0, unsigned long id1, unsigned long size0, unsigned long size1) {
  g_item.global_id[0] = id0;
  g_item.global_id[1] = id1;
  g_item.global_size[0] = size0;
  g_item.global_size[1] = size1;
}

int fiber_lane() { return g_group ? g_group->cur : 0; }

void fiber_yield() {
  Group *g = g_group;
  if (_setjmp(g->lane[g->cur].ctx) == 0) _longjmp(g->sched, 1);
}

void run_workgroup(void (*body)(void *), void *arg, int lanes) {
  Group *g = new Group();
  g->nlanes = lanes;
  g->body = body;
  g->arg = arg;
  Group *saved = g_group;
  g_group = g;
  for (int i = 0; i < lanes; i++) {
    Lane &l = g->lane[i];
    l.stack = (char *)malloc(kStack);
    l.done = false;
    getcontext(&l.boot);
    l.boot.uc_stack.ss_sp = l.stack;
    l.boot.uc_stack.ss_size = kStack;
    l.boot.uc_link = nullptr;
    makecontext(&l.boot, (void (*)())trampoline, 0);
    g->cur = i;
    if (_setjmp(g->sched) == 0) swapcontext(&g->sched_uc, &l.boot);
  }
  /* round robin: one pass over the lanes is one barrier phase */
  for (;;) {
    int alive = 0;
    for (int i = 0; i < lanes; i++) {
      if (g->lane[i].done) continue;
      g->cur = i;
      if (_setjmp(g->sched) == 0) _longjmp(g->lane[i].ctx, 1);
      alive += !g->lane[i].done;
    }
    if (!alive) break;
  }
  for (int i = 0; i < lanes; i++) free(g->lane[i].stack);
  g_group = saved;
  delete g;
}

}  // namespace refshim
