// Shared by the five command lines: the reference's timer (core/time.hpp:22-26)
// and its "active(i)>=n" lines, rebuilt from the per-call trace.
#ifndef GEMINI_GB300_TOOLKIT_COMMON_HPP
#define GEMINI_GB300_TOOLKIT_COMMON_HPP

#include <stdio.h>
#include <stdlib.h>
#include <sys/time.h>

#include "gemini/graph.hpp"

inline double get_time() {
  struct timeval tv;
  gettimeofday(&tv, NULL);
  return tv.tv_sec + (tv.tv_usec / 1e6);
}

// The reference prints, at the top of iteration i, the count its previous
// process_edges call activated (first: `first`) for calls [0, calls).
inline void print_active(const TraceBuffers &tb, int calls, unsigned long long first) {
  unsigned long long active = first;
  for (int i = 0; i < calls; i++) {
    printf("active(%d)>=%llu\n", i, active);
    active = tb.activated[i];
  }
}

template <typename F>
int run_main(F body) {
  try {
    body();
  } catch (const gemini::Error &e) {
    fprintf(stderr, "%s\n", e.what());
    return 1;
  }
  return 0;
}

#endif
