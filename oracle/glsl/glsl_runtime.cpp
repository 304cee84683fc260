// TEST INFRASTRUCTURE ONLY — the dispatch loop of the host GLSL environment (glsl.hpp).
//
// A dispatch runs its workgroups one after the other.  The first invocation of the dispatch runs
// on a fiber: if it finishes without reaching barrier(), the shader takes no workgroup-wide step
// on this dispatch (barriers sit in uniform control flow), and every other invocation runs to
// completion in turn.  If it reaches a barrier, every workgroup of the dispatch runs its 128
// invocations as fibers, each resumed in turn until the next barrier, so that all of them
// reach a barrier before any passes it.
#include <ucontext.h>

#include <cstdio>
#include <cstdlib>
#include <vector>

#include "glsl.hpp"

namespace glsl {

Invocation* current = nullptr;

namespace {

constexpr int kLocal = 128;
constexpr size_t kStack = 256 * 1024;

struct Fiber {
  ucontext_t ctx;
  Invocation inv;
  bool done = false;
  bool waiting = false;
  std::vector<char> stack;
};

ucontext_t g_scheduler;
Fiber* g_running = nullptr;  // the fiber being resumed, null when running directly
void (*g_body)() = nullptr;
std::vector<Fiber> g_fibers;

void run_fiber() {
  g_body();
  g_running->done = true;
  // returning resumes uc_link (the scheduler)
}

void start(Fiber& f, const Invocation& inv) {
  f.inv = inv;
  f.done = false;
  f.waiting = false;
  if (f.stack.empty()) f.stack.resize(kStack);
  getcontext(&f.ctx);
  f.ctx.uc_stack.ss_sp = f.stack.data();
  f.ctx.uc_stack.ss_size = f.stack.size();
  f.ctx.uc_link = &g_scheduler;
  makecontext(&f.ctx, run_fiber, 0);
}

// Resumes f until it finishes or reaches a barrier.
void resume(Fiber& f) {
  g_running = &f;
  current = &f.inv;
  f.waiting = false;
  swapcontext(&g_scheduler, &f.ctx);
  g_running = nullptr;
}

Invocation make(uvec3 groups, uint gx, uint gy, uint lid) {
  Invocation inv;
  inv.groups = groups;
  inv.group = uvec3(gx, gy, 0u);
  inv.local = uvec3(lid, 0u, 0u);
  inv.global = uvec3(gx * kLocal + lid, gy, 0u);
  return inv;
}

// All 128 invocations of one workgroup as fibers; fiber 0 may already have started.
void run_group_fibers(uvec3 groups, uint gx, uint gy, bool first_started) {
  for (int k = 0; k < kLocal; k++)
    if (!(k == 0 && first_started)) start(g_fibers[k], make(groups, gx, gy, (uint)k));
  // a first fiber that already waits at its first barrier stays there until the others reach it
  if (first_started)
    for (int k = 1; k < kLocal; k++) resume(g_fibers[k]);
  int live = 0;
  for (int k = 0; k < kLocal; k++) live += g_fibers[k].done ? 0 : 1;
  while (live > 0) {
    for (int k = 0; k < kLocal; k++) {
      Fiber& f = g_fibers[k];
      if (f.done) continue;
      resume(f);
      if (f.done) live--;
    }
  }
}

}  // namespace

void barrier() {
  if (!g_running) {
    std::fprintf(stderr, "glsl: barrier() outside a fiber (non-uniform barrier in a dispatch)\n");
    std::abort();
  }
  Fiber* f = g_running;
  f->waiting = true;
  swapcontext(&f->ctx, &g_scheduler);
}

void dispatch(void (*body)(), uvec3 groups) {
  if (g_fibers.size() < (size_t)kLocal) g_fibers.resize(kLocal);
  g_body = body;
  if (groups.x == 0 || groups.y == 0) return;
  // probe: invocation 0 of workgroup 0 on a fiber
  start(g_fibers[0], make(groups, 0, 0, 0));
  resume(g_fibers[0]);
  const bool cooperative = !g_fibers[0].done;
  for (uint gy = 0; gy < groups.y; gy++)
    for (uint gx = 0; gx < groups.x; gx++) {
      const bool first = gx == 0 && gy == 0;
      if (cooperative) {
        run_group_fibers(groups, gx, gy, first);
        continue;
      }
      for (uint lid = first ? 1u : 0u; lid < (uint)kLocal; lid++) {
        Invocation inv = make(groups, gx, gy, lid);
        current = &inv;
        body();
      }
    }
  current = nullptr;
}

}  // namespace glsl
