// Host check of the pool's free-extent bookkeeping (anuga_core_gb300/csrc/
// free_runs.h) against a plain owner array scanned the way the pool once did:
// random allocations (first fit: the lowest free run that fits) and releases
// of scenario-sized extents; after every operation the two agree on where an
// extent goes, the largest free run and one past the last used unit.
//   check_free_runs [operations]
#include <cstdio>
#include <cstdlib>
#include <random>
#include <vector>
#include "../../anuga_core_gb300/csrc/free_runs.h"

static long long first_fit(const std::vector<int>& own, long long len) {
  long long run = 0;
  for (long long i = 0; i < (long long)own.size(); i++) {
    run = own[i] < 0 ? run + 1 : 0;
    if (run == len) return i - len + 1;
  }
  return -1;
}
static long long largest(const std::vector<int>& own) {
  long long run = 0, m = 0;
  for (int o : own) { run = o < 0 ? run + 1 : 0; m = std::max(m, run); }
  return m;
}
static long long used_end(const std::vector<int>& own) {
  long long e = 0;
  for (long long i = 0; i < (long long)own.size(); i++) if (own[i] >= 0) e = i + 1;
  return e;
}

int main(int argc, char** argv) {
  const long long ops = argc > 1 ? std::atoll(argv[1]) : 20000;
  std::mt19937_64 rng(7);
  long long bad = 0;
  for (int trial = 0; trial < 4; trial++) {
    const long long n = 200 + 300 * trial;
    std::vector<int> own(n, -1);
    agx::FreeRuns fr;
    fr.init(n);
    std::vector<std::pair<long long, long long>> live;        // (start, len)
    for (long long op = 0; op < ops; op++) {
      const bool add = live.empty() || (rng() % 100) < 55;
      if (add) {
        const long long len = 1 + (long long)(rng() % (1 + n / (4 + rng() % 12)));
        const long long a = first_fit(own, len), b = fr.find(len);
        if (a != b) bad++;
        if (a >= 0) {
          for (long long i = a; i < a + len; i++) own[i] = 1;
          fr.take(a, len);
          live.push_back({a, len});
        }
      } else {
        const size_t k = rng() % live.size();
        const auto e = live[k];
        live.erase(live.begin() + k);
        for (long long i = e.first; i < e.first + e.second; i++) own[i] = -1;
        fr.give(e.first, e.second);
      }
      if (largest(own) != fr.largest() || used_end(own) != fr.used_end()) bad++;
    }
  }
  std::printf("mismatches %lld\n", bad);
  return bad ? 1 : 0;
}
