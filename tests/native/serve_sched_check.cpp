// Checks of the request server's host bookkeeping (serve_sched.h): slot
// arena against a bitmap model under random alloc/release sequences, the
// admission order with backfilling and its bypass bound, and percentiles.
#include <cstdio>
#include <cstdlib>
#include <random>

#include "serve_sched.h"

using namespace gbrkc::serve;

static int failures = 0;
#define CHECK(c)                                                   \
  do {                                                             \
    if (!(c)) {                                                    \
      std::printf("FAIL %s:%d: %s\n", __FILE__, __LINE__, #c);     \
      failures++;                                                  \
    }                                                              \
  } while (0)

static void arena_basics() {
  SlotArena a(10);
  std::vector<Run> r1, r2, r3, r4;
  CHECK(a.alloc(4, r1) && r1.size() == 1 && r1[0] == Run(0, 4));
  CHECK(a.alloc(3, r2) && r2[0] == Run(4, 3));
  CHECK(a.alloc(3, r3) && r3[0] == Run(7, 3));
  CHECK(a.free_slots() == 0 && !a.alloc(1, r4) && r4.empty());
  a.release(r1);
  a.release(r3);
  CHECK(a.free_slots() == 7 && a.gaps() == 2);
  // no gap of 5: two runs in address order
  CHECK(a.alloc(5, r4) && r4.size() == 2 && r4[0] == Run(0, 4) && r4[1] == Run(7, 1));
  a.release(r4);
  a.release(r2);
  CHECK(a.free_slots() == 10 && a.gaps() == 1);
  std::vector<Run> r5;
  CHECK(!a.alloc(11, r5) && a.free_slots() == 10);
  CHECK(!a.alloc(0, r5));
}

static void arena_random() {
  std::mt19937 rng(12345);
  const int N = 257;
  SlotArena a(N);
  std::vector<int> used(N, -1);
  std::vector<std::vector<Run>> live;
  for (int step = 0; step < 20000; step++) {
    if (!live.empty() && (rng() % 3 == 0 || a.free_slots() == 0)) {
      const size_t k = rng() % live.size();
      for (const Run &r : live[k])
        for (int i = r.first; i < r.first + r.second; i++) {
          CHECK(used[i] >= 0);
          used[i] = -1;
        }
      a.release(live[k]);
      live.erase(live.begin() + k);
    } else {
      const int n = 1 + rng() % 40;
      std::vector<Run> runs;
      const int before = a.free_slots();
      const bool ok = a.alloc(n, runs);
      CHECK(ok == (n <= before));
      if (!ok) continue;
      int got = 0;
      for (const Run &r : runs) {
        CHECK(r.second > 0 && r.first >= 0 && r.first + r.second <= N);
        for (int i = r.first; i < r.first + r.second; i++) {
          CHECK(used[i] < 0);
          used[i] = step;
        }
        got += r.second;
      }
      CHECK(got == n && a.free_slots() == before - n);
      live.push_back(runs);
    }
    int fr = 0;
    for (int u : used) fr += (u < 0);
    CHECK(fr == a.free_slots());
  }
  for (auto &r : live) a.release(r);
  CHECK(a.free_slots() == N && a.gaps() == 1);
}

static void admission() {
  // sizes of requests 0..4 against 10 free units
  std::vector<int> size = {6, 8, 3, 2, 5};
  int free_units = 10;
  Admission q(2);
  for (int i = 0; i < 5; i++) q.push(i);
  auto fits = [&](int r) {
    if (size[r] > free_units) return false;
    free_units -= size[r];
    return true;
  };
  std::vector<int> a = q.admit(fits);  // 0 (6), head 1 (8) does not fit; backfill 2 (3)
  CHECK(a.size() == 2 && a[0] == 0 && a[1] == 2 && free_units == 1);
  free_units += 6;  // request 0 done: 7 free; head 1 still does not fit; 3 (2) and 4 (5) do
  a = q.admit(fits);
  CHECK(a.size() == 2 && a[0] == 3 && a[1] == 4 && free_units == 0 && q.size() == 1);
  // the head has now been passed over twice: nothing overtakes it any more
  q.push(5);
  size.push_back(1);
  free_units = 1;
  a = q.admit(fits);
  CHECK(a.empty() && q.size() == 2);
  free_units = 9;
  a = q.admit(fits);
  CHECK(a.size() == 2 && a[0] == 1 && a[1] == 5 && q.empty());
  Admission r;
  r.push(7);
  r.push(8);
  CHECK(r.remove(7) && !r.remove(7) && r.size() == 1);
}

static void percentiles() {
  std::vector<double> v;
  for (int i = 1; i <= 100; i++) v.push_back(101 - i);
  CHECK(percentile(v, 50) == 50.0 && percentile(v, 99) == 99.0 && percentile(v, 100) == 100.0);
  CHECK(percentile(v, 0) == 1.0);
  CHECK(percentile({}, 50) == 0.0);
  CHECK(percentile({3.0}, 99) == 3.0);
}

int main() {
  arena_basics();
  arena_random();
  admission();
  percentiles();
  if (failures) return 1;
  std::printf("OK\n");
  return 0;
}
