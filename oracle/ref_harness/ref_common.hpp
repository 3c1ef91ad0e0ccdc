/* Shared helpers for the reference-program harnesses (oracle/_ref/*).
 * Test infrastructure: these mains drive the reference's own CPU functions,
 * compiled from its sources in place, and dump per-vertex results in binary. */
#pragma once
#include <chrono>
#include <climits>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iomanip>
#include <iostream>
#include <map>
#include <string>
#include <vector>
#include <ctime>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

static inline uint64_t og_ref_read_vertex_count(const char *path) {
  uint64_t v = 0;
  FILE *f = fopen(path, "rb");
  if (!f || fread(&v, 8, 1, f) != 1) {
    fprintf(stderr, "cannot read %s\n", path);
    exit(2);
  }
  fclose(f);
  return v;
}

static inline void og_ref_write(const char *path, const void *p, size_t n) {
  FILE *f = fopen(path, "ab");
  if (!f || fwrite(p, 1, n, f) != n) {
    fprintf(stderr, "cannot write %s\n", path);
    exit(2);
  }
  fclose(f);
}

static inline double og_ref_now_ms() {
  return std::chrono::duration<double, std::milli>(
             std::chrono::steady_clock::now().time_since_epoch())
      .count();
}
