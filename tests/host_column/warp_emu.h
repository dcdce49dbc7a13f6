// TEST INFRASTRUCTURE -- not part of the product and never loaded by it.
//
// A 32-lane warp on one host thread, for running the product's warp-cooperative
// device code on the CPU.  Each lane is a fiber (ucontext) running the same function;
// a lane runs until its next warp collective (__syncwarp, a shuffle, a ballot), which
// is a barrier: when every lane has arrived the collective's results are formed and
// the lanes resume, each round in a fresh seeded random order.  Memory written by
// one lane between two collectives is therefore seen by the others in an order that
// changes from round to round, so device code that reads another lane's writes
// without a barrier in between gives results that depend on the seed.
//
// Requires every lane to call the same collectives in the same order (full-mask,
// convergent use, which is how the device code uses them); run() reports a mismatch.

#pragma once

#include <ucontext.h>

#include <algorithm>
#include <cstdint>
#include <functional>
#include <random>
#include <vector>

namespace warp_emu {

enum Kind { kSync = 1, kShfl = 2, kShflUp = 3, kBallot = 4, kShflXor = 5, kMatch = 6 };

struct Warp {
  ucontext_t sched;
  ucontext_t ctx[32];
  std::vector<char> stack[32];
  void* schedJmp[5];    // __builtin_setjmp buffers: switching lanes this way keeps the
  void* laneJmp[32][5];  // signal mask alone (swapcontext makes a system call each time)
  bool started[32];
  bool finished[32];
  int kind[32];
  uint32_t value[32];
  int arg[32];
  uint32_t result[32];
  const std::function<void(int)>* body;
  int lane;
};

inline thread_local Warp* g_warp = nullptr;

// (a function may not both __builtin_setjmp and __builtin_longjmp: each jump has its own)
__attribute__((noinline)) inline void jumpScheduler(Warp* w) { __builtin_longjmp(w->schedJmp, 1); }

__attribute__((noinline)) inline void jumpLane(Warp* w, int lane) {
  if (w->started[lane]) __builtin_longjmp(w->laneJmp[lane], 1);
  w->started[lane] = true;
  setcontext(&w->ctx[lane]);  // first entry onto the fiber's own stack
}

__attribute__((noinline)) inline void toScheduler(Warp* w, int lane) {
  if (__builtin_setjmp(w->laneJmp[lane]) == 0) jumpScheduler(w);
}

__attribute__((noinline)) inline void toLane(Warp* w, int lane) {
  if (__builtin_setjmp(w->schedJmp) == 0) jumpLane(w, lane);
}

inline void trampoline() {
  Warp* w = g_warp;
  const int lane = w->lane;
  (*w->body)(lane);
  w->finished[lane] = true;
  jumpScheduler(w);
}

inline uint32_t collective(int kind, uint32_t v, int arg) {
  Warp* w = g_warp;
  const int lane = w->lane;
  w->kind[lane] = kind;
  w->value[lane] = v;
  w->arg[lane] = arg;
  toScheduler(w, lane);
  return w->result[lane];
}

// Runs body(lane) for lanes 0..31.  Returns false when the lanes' collectives did not
// match (different kinds at one barrier, or some lanes finished while others wait).
inline bool run(const std::function<void(int)>& body, uint64_t seed) {
  Warp w;
  Warp* saved = g_warp;
  g_warp = &w;
  w.body = &body;
  for (int l = 0; l < 32; ++l) {
    w.stack[l].resize(1 << 18);
    getcontext(&w.ctx[l]);
    w.ctx[l].uc_stack.ss_sp = w.stack[l].data();
    w.ctx[l].uc_stack.ss_size = w.stack[l].size();
    w.ctx[l].uc_link = &w.sched;
    makecontext(&w.ctx[l], trampoline, 0);
    w.started[l] = false;
    w.finished[l] = false;
  }
  std::mt19937_64 rng(seed);
  int order[32];
  for (int l = 0; l < 32; ++l) order[l] = l;
  bool ok = true;
  for (;;) {
    std::shuffle(order, order + 32, rng);
    for (int i = 0; i < 32; ++i) {
      const int l = order[i];
      if (w.finished[l]) continue;
      w.lane = l;
      toLane(&w, l);
    }
    int done = 0;
    for (int l = 0; l < 32; ++l) done += w.finished[l] ? 1 : 0;
    if (done == 32) break;
    if (done != 0) {
      ok = false;
      break;
    }
    const int kind = w.kind[0];
    for (int l = 1; l < 32; ++l)
      if (w.kind[l] != kind) ok = false;
    if (!ok) break;
    uint32_t ballot = 0;
    for (int l = 0; l < 32; ++l)
      if (w.value[l]) ballot |= 1u << l;
    for (int l = 0; l < 32; ++l) {
      switch (kind) {
        case kShfl: w.result[l] = w.value[w.arg[l] & 31]; break;
        case kShflUp: w.result[l] = l - w.arg[l] >= 0 ? w.value[l - w.arg[l]] : w.value[l]; break;
        case kBallot: w.result[l] = ballot; break;
        case kShflXor: w.result[l] = w.value[(l ^ w.arg[l]) & 31]; break;
        case kMatch: {
          uint32_t m = 0;
          for (int o = 0; o < 32; ++o)
            if (w.value[o] == w.value[l]) m |= 1u << o;
          w.result[l] = m;
          break;
        }
        default: w.result[l] = 0; break;
      }
    }
  }
  g_warp = saved;
  return ok;
}

}  // namespace warp_emu
